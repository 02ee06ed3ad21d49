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

# The "Mode6Index2 fast" variant (oracle/ref_m6i2_only.cpp): the mode files'
# own fast passes renamed away, empty ones linked in their place; the
# preset is the default one (Mode6Index2 runs only with kDenoise or
# kDenoiseStep non-zero, src/Bc7Core.cpp:1548).
D=1; S=9
LIB="$OUT/libnebc7_ref_d${D}s${S}_m6i2.so"
OBJ="$OUT/obj_d${D}s${S}_m6i2"
mkdir -p "$OBJ"
pids=""
for f in $FILES; do
  EXTRA=""
  case "$f" in
    Bc7CoreMode6Index2.cpp) ;;
    Bc7CoreMode*.cpp) EXTRA="-DCompressBlockFast=CompressBlockFastOff" ;;
  esac
  g++ -O2 -std=c++17 -mavx2 -mfma -mbmi -mbmi2 -mlzcnt -mpopcnt -ffp-contract=off \
    -fPIC -w -DOPTION_LIBRARY -DNEBC7_REF_DENOISE=$D -DNEBC7_REF_DENOISE_STEP=$S $EXTRA \
    -include "$HERE/ref_shim.h" -I"$SRC" -c "$SRC/$f" -o "$OBJ/${f%.cpp}.o" &
  pids="$pids $!"
done
for extra in ref_harness ref_m6i2_only; do
  g++ -O2 -std=c++17 -mavx2 -mfma -mbmi -mbmi2 -mlzcnt -mpopcnt -ffp-contract=off \
    -fPIC -w -DOPTION_LIBRARY -DNEBC7_REF_DENOISE=$D -DNEBC7_REF_DENOISE_STEP=$S \
    -include "$HERE/ref_shim.h" -I"$SRC" -c "$HERE/$extra.cpp" -o "$OBJ/$extra.o" &
  pids="$pids $!"
done
for p in $pids; do wait $p; done
g++ -shared -o "$LIB" "$OBJ"/*.o -lpthread
echo "built $LIB"

# The command-line build (oracle/ref_cli_shim.h, ref_cli_harness.cpp): every
# source with the reference's own configuration (src/Bc7Mode.h) and without
# OPTION_LIBRARY, for the CLI's /map and /bad outputs and its real job pool.
LIB="$OUT/libnebc7_ref_cli.so"
OBJ="$OUT/obj_cli"
mkdir -p "$OBJ"
pids=""
# -fno-semantic-interposition: gcc refuses the reference's always_inline on
# functions it may interpose under -fPIC (src/pch.h:34-37 omits `inline`)
for f in $FILES Worker.cpp; do
  g++ -O2 -std=c++17 -mavx2 -mfma -mbmi -mbmi2 -mlzcnt -mpopcnt -ffp-contract=off \
    -fPIC -fno-semantic-interposition -w -include "$HERE/ref_cli_shim.h" -I"$SRC" -c "$SRC/$f" -o "$OBJ/${f%.cpp}.o" &
  pids="$pids $!"
done
g++ -O2 -std=c++17 -mavx2 -mfma -mbmi -mbmi2 -mlzcnt -mpopcnt -ffp-contract=off \
  -fPIC -fno-semantic-interposition -w -include "$HERE/ref_cli_shim.h" -I"$SRC" -c "$HERE/ref_cli_harness.cpp" -o "$OBJ/ref_cli_harness.o" &
pids="$pids $!"
for p in $pids; do wait $p; done
# header functions marked always_inline without `inline` (src/Bc7Core.h:123
# GetArea) are emitted by every file that includes them: identical copies
g++ -shared -Wl,-z,muldefs -o "$LIB" "$OBJ"/*.o -lpthread
echo "built $LIB"
