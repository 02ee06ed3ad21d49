#!/bin/sh
# Builds the reference encoder from its own sources as the CPU oracle
# (test infrastructure only).  Output goes to oracle/_ref/ (git-ignored).
# The sources are read where they lie; nothing is copied into this repository.
#
#   usage: oracle/build_ref.sh [reference_src_dir]
#
# Without an argument the sources are taken from $NEBC7_REFERENCE_SRC, else
# from a checkout named `reference` beside this repository.
#
# One shared library per (kDenoise, kDenoiseStep) preset, because the
# reference fixes the preset at compile time (src/Bc7Mode.h:10-13).
# -ffp-contract=off keeps the double-precision SSIM tie-break
# (src/Bc7Core.cpp:1341-1428) unfused, as the reference's MSVC build computes it.
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
SRC=${1:-${NEBC7_REFERENCE_SRC:-$HERE/../../reference/src}}
OUT="$HERE/_ref"
if [ ! -d "$SRC" ]; then
  echo "reference sources not found at $SRC; skipping" >&2
  exit 0
fi
case "$(uname -m)" in
  x86_64|amd64) ;;
  *) echo "reference build needs x86-64 SIMD; skipping on $(uname -m)" >&2; exit 0 ;;
esac
mkdir -p "$OUT"
FILES="Bc7Core.cpp Bc7Tables.cpp Metrics.cpp Bc7Compress.cpp \
  Bc7CoreMode0.cpp Bc7CoreMode1.cpp Bc7CoreMode2.cpp Bc7CoreMode3.cpp \
  Bc7CoreMode4.cpp Bc7CoreMode5.cpp Bc7CoreMode6.cpp Bc7CoreMode6Index2.cpp Bc7CoreMode7.cpp"
for preset in "1 9" "0 0" "1 0" "0 9"; do
  set -- $preset
  D=$1; S=$2
  LIB="$OUT/libnebc7_ref_d${D}s${S}.so"
  OBJ="$OUT/obj_d${D}s${S}"
  mkdir -p "$OBJ"
  pids=""
  for f in $FILES; do
    g++ -O2 -std=c++17 -mavx2 -mfma -mbmi -mbmi2 -mlzcnt -mpopcnt -ffp-contract=off \
      -fPIC -w -DOPTION_LIBRARY -DNEBC7_REF_DENOISE=$D -DNEBC7_REF_DENOISE_STEP=$S \
      -include "$HERE/ref_shim.h" -I"$SRC" -c "$SRC/$f" -o "$OBJ/${f%.cpp}.o" &
    pids="$pids $!"
  done
  g++ -O2 -std=c++17 -mavx2 -mfma -mbmi -mbmi2 -mlzcnt -mpopcnt -ffp-contract=off \
    -fPIC -w -DOPTION_LIBRARY -DNEBC7_REF_DENOISE=$D -DNEBC7_REF_DENOISE_STEP=$S \
    -include "$HERE/ref_shim.h" -I"$SRC" -c "$HERE/ref_harness.cpp" -o "$OBJ/ref_harness.o" &
  pids="$pids $!"
  for p in $pids; do wait $p; done
  g++ -shared -o "$LIB" "$OBJ"/*.o -lpthread
  echo "built $LIB"
done
